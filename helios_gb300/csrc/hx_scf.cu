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
#include "hx_common.cuh"
#include "hx_plan.h"

namespace {
constexpr int NT = 512;

__device__ double block_reduce(double v, double *sh, bool is_max)
{
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = is_max ? fmax(v, w) : v + w;
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : (is_max ? 0.0 : 0.0);
        for (int o = 16; o > 0; o >>= 1) {
            double w = __shfl_xor_sync(0xffffffffu, v, o);
            v = is_max ? fmax(v, w) : v + w;
        }
        if (lane == 0) sh[32] = v;
    }
    __syncthreads();
    double r = sh[32];
    __syncthreads();
    return r;
}

// C = op(A) op(B) for N x N row-major matrices (ta/tb: use the transpose).
__device__ void mm(double *C, const double *A, const double *B, int n, bool ta, bool tb, int kmax)
{
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int i = e / n, j = e % n;
        double s = 0.0;
        for (int k = 0; k < kmax; ++k) {
            double a = ta ? A[k * n + i] : A[i * n + k];
            double b = tb ? B[j * n + k] : B[k * n + j];
            s = fma(a, b, s);
        }
        C[e] = s;
    }
    __syncthreads();
}

// F = core - G o D + 2 diag(G diag D)
__device__ void fock(double *F, const double *core, const double *G, const double *D, int n)
{
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int i = e / n, j = e % n;
        double f = core[e] - G[e] * D[e];
        if (i == j) {
            double s = 0.0;
            for (int l = 0; l < n; ++l) s += G[i * n + l] * D[l * n + l];
            f += 2.0 * s;
        }
        F[e] = f;
    }
    __syncthreads();
}

// D = sum_{i<nocc} V[:,i] V[:,i]^T
__device__ void density(double *D, const double *V, int n, int nocc)
{
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int mu = e / n, nu = e % n;
        double s = 0.0;
        for (int i = 0; i < nocc; ++i) s = fma(V[mu * n + i], V[nu * n + i], s);
        D[e] = s;
    }
    __syncthreads();
}

// Jacobi eigen-decomposition of symmetric A (n x n, destroyed: its diagonal
// ends as the eigenvalues); rotations accumulate into V. W is n x n scratch.
// Afterwards V's columns and E are sorted ascending.
__device__ int jacobi(double *A, double *V, double *E, double *W, int n, double *sh,
                      int *pp, int *pq, double *pc, double *ps)
{
    const int np = n + (n & 1);
    int sweeps = 0;
    for (; sweeps < 40; ++sweeps) {
        double off = 0.0, tot = 0.0;
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            double a = A[e] * A[e];
            tot += a;
            if (e / n != e % n) off += a;
        }
        off = block_reduce(off, sh, false);
        tot = block_reduce(tot, sh, false);
        if (off <= 1e-30 * tot || off < 1e-300) break;
        for (int r = 0; r < np - 1; ++r) {
            for (int k = threadIdx.x; k < np / 2; k += blockDim.x) {
                int x = k, y = np - 1 - k;
                int p = (x == 0) ? 0 : 1 + (x - 1 + r) % (np - 1);
                int q = 1 + (y - 1 + r) % (np - 1);
                if (p > q) { int t = p; p = q; q = t; }
                double c = 1.0, s = 0.0;
                if (q < n) {
                    double apq = A[p * n + q];
                    if (fabs(apq) > 1e-300) {
                        double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                        double t;
                        if (fabs(theta) > 1e150) t = 0.5 / theta;
                        else t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0);
                        s = t * c;
                    }
                } else {
                    p = -1;   // bye for odd n
                }
                pp[k] = p; pq[k] = q; pc[k] = c; ps[k] = s;
            }
            __syncthreads();
            // columns of A and V: X <- X J
            for (int e = threadIdx.x; e < (np / 2) * n; e += blockDim.x) {
                int k = e / n, row = e % n, p = pp[k], q = pq[k];
                if (p < 0 || ps[k] == 0.0) continue;
                double c = pc[k], s = ps[k];
                double akp = A[row * n + p], akq = A[row * n + q];
                A[row * n + p] = c * akp - s * akq;
                A[row * n + q] = s * akp + c * akq;
                double vkp = V[row * n + p], vkq = V[row * n + q];
                V[row * n + p] = c * vkp - s * vkq;
                V[row * n + q] = s * vkp + c * vkq;
            }
            __syncthreads();
            // rows of A: A <- J^T A
            for (int e = threadIdx.x; e < (np / 2) * n; e += blockDim.x) {
                int k = e / n, col = e % n, p = pp[k], q = pq[k];
                if (p < 0 || ps[k] == 0.0) continue;
                double c = pc[k], s = ps[k];
                double apk = A[p * n + col], aqk = A[q * n + col];
                A[p * n + col] = c * apk - s * aqk;
                A[q * n + col] = s * apk + c * aqk;
            }
            __syncthreads();
        }
    }
    // sort ascending: rank each eigenvalue, permute V's columns through W
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
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
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) V[e] = W[e];
    __syncthreads();
    return sweeps;
}

__global__ void __launch_bounds__(NT) scf_kernel(const ScfMol *__restrict__ mols, ScfParams prm)
{
    __shared__ double sh[40];
    __shared__ int pp[HX_MAX_MOL_N / 2], pq[HX_MAX_MOL_N / 2];
    __shared__ double pc[HX_MAX_MOL_N / 2], ps[HX_MAX_MOL_N / 2];
    const ScfMol m = mols[blockIdx.x];
    const int n = m.N, no = m.nocc, nn = n * n;
    double *F = m.F, *D = m.D, *V = m.V, *A = m.A, *W1 = m.W1, *W2 = m.W2;

    // guess
    if (m.D0) {
        for (int e = threadIdx.x; e < nn; e += blockDim.x) D[e] = m.D0[e];
        for (int e = threadIdx.x; e < nn; e += blockDim.x) V[e] = m.V0 ? m.V0[e] : (e / n == e % n);
        __syncthreads();
    } else {
        for (int e = threadIdx.x; e < nn; e += blockDim.x) {
            A[e] = m.huckel[e];
            V[e] = (e / n == e % n) ? 1.0 : 0.0;
        }
        __syncthreads();
        jacobi(A, V, m.E, W1, n, sh, pp, pq, pc, ps);
        density(D, V, n, no);
    }
    fock(F, m.core, m.G, D, n);

    int iteration = 0, successful = 1, status = 0;
    double current = 0.0;
    for (;;) {
        ++iteration;
        // W1 = F R, R = 2D - 1
        for (int e = threadIdx.x; e < nn; e += blockDim.x) W2[e] = 2.0 * D[e] - (e / n == e % n);
        __syncthreads();
        mm(W1, F, W2, n, false, false, n);
        // A = W1 - W1^T  (F R - R F, both symmetric)
        for (int e = threadIdx.x; e < nn; e += blockDim.x) A[e] = W1[e] - W1[(e % n) * n + e / n];
        __syncthreads();
        mm(W1, A, W2, n, false, false, n);           // Fmin
        double acc = 0.0;
        for (int e = threadIdx.x; e < nn; e += blockDim.x) acc = fmax(acc, fabs(W1[e]));
        acc = block_reduce(acc, sh, true);
        for (int e = threadIdx.x; e < nn; e += blockDim.x) D[e] -= prm.step * W1[e];
        __syncthreads();
        fock(F, m.core, m.G, D, n);
        // diagonalise F in the current basis: A = V^T F V
        mm(W1, F, V, n, false, false, n);
        mm(A, V, W1, n, true, false, n);
        jacobi(A, V, m.E, W1, n, sh, pp, pq, pc, ps);
        density(D, V, n, no);
        fock(F, m.core, m.G, D, n);

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
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        eel += D[e] * (m.core[e] + F[e]);
        if (e / n < e % n) enuc += m.G[e];
    }
    eel = block_reduce(eel, sh, false);
    enuc = block_reduce(enuc, sh, false);
    if (threadIdx.x == 0) {
        m.out[0] = eel + enuc;
        m.out[1] = eel;
        m.out[2] = enuc;
        m.out[3] = current;
        m.status[0] = status;
        m.status[1] = iteration;
    }
}

// MO Fock (prepareFock('spatial'), mod_cc.f90:2336-2396): Fmo = V^T F V.
__global__ void __launch_bounds__(NT) mo_fock_kernel(const ScfMol *__restrict__ mols)
{
    const ScfMol m = mols[blockIdx.x];
    mm(m.W1, m.F, m.V, m.N, false, false, m.N);
    mm(m.Fmo, m.V, m.W1, m.N, true, false, m.N);
}
}  // namespace

cudaError_t hx_scf_launch(const ScfMol *d_mols, int nmol, const ScfParams &p, cudaStream_t s)
{
    scf_kernel<<<nmol, NT, 0, s>>>(d_mols, p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    mo_fock_kernel<<<nmol, NT, 0, s>>>(d_mols);
    return cudaGetLastError();
}
