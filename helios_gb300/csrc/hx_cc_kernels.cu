// Elementwise, reduction and DIIS kernels of the CCSD iteration (FP64, HBM bound).
//
// All kernels are grouped over the molecules of a batch: blockIdx.y selects
// the molecule, blockIdx.x strides over its elements, and molecules whose
// `active` flag is 0 return at once. Reductions are two-pass (fixed per-block
// partials, then an ordered sum), so repeated runs are bitwise identical.
#include "hx_common.cuh"
#include "hx_plan.h"
#include "hx_kernels.h"

namespace {
constexpr int NT = 256;

__device__ __forceinline__ bool skip(const int *active) { return active && !active[blockIdx.y]; }

#define GRID_LOOP(i, n) for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
                             i += (long long)gridDim.x * blockDim.x)

__device__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ double warp_max(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
// block-wide reduction (sum or max) of blockDim.x == NT threads
__device__ double block_red(double v, bool mx)
{
    __shared__ double sh[NT / 32];
    v = mx ? warp_max(v) : warp_sum(v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    v = (threadIdx.x < NT / 32) ? sh[threadIdx.x] : 0.0;
    if (w == 0) v = mx ? warp_max(v) : warp_sum(v);
    return v;   // valid in thread 0
}

// ---------------------------------------------------------------- dressing
// X = [Co | Cv], Y = [Co | Cv]; the t1 corrections are added by GEMMs.
__global__ void k_dress_init(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const long long nn = (long long)m.N * m.N;
    GRID_LOOP(e, nn) { m.X[e] = m.Cmo[e]; m.Y[e] = m.Cmo[e]; }
}

// H2 = h - G o Pm + 2 diag(G diag Pm), Pm = Yo Xo^T (dressed half density)
__global__ void k_dress_fock(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int n = m.N;
    GRID_LOOP(e, (long long)n * n) {
        int i = (int)(e / n), j = (int)(e % n);
        double f = m.h[e] - m.G[e] * m.Pm[e];
        if (i == j) {
            double s = 0.0;
            for (int l = 0; l < n; ++l) s += m.G[i * n + l] * m.Pm[l * n + l];
            f += 2.0 * s;
        }
        m.H2[e] = f;
    }
}

// ZDO pair products of the dressed factors.
__global__ void k_zdo_products(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int n = m.N, o = m.o, v = m.v;
    const long long nia = (long long)n * o * v, noo = (long long)n * o * o, nvv = (long long)n * v * v;
    GRID_LOOP(e, nia + noo + nvv) {
        if (e < nia) {
            int mu = (int)(e / (o * v)), r = (int)(e % (o * v)), i = r / v, a = r % v;
            m.Bia[e] = m.X[mu * n + o + a] * m.Y[mu * n + i];
        } else if (e < nia + noo) {
            long long f = e - nia;
            int mu = (int)(f / (o * o)), r = (int)(f % (o * o)), k = r / o, i = r % o;
            m.Boo[f] = m.X[mu * n + k] * m.Y[mu * n + i];
        } else {
            long long f = e - nia - noo;
            int mu = (int)(f / (v * v)), r = (int)(f % (v * v)), a = r / v, c = r % v;
            m.Bvv[f] = m.X[mu * n + o + a] * m.Y[mu * n + o + c];
        }
    }
}

// u[i][a][j][b] = 2 t[i][a][j][b] - t[i][b][j][a]
__global__ void k_make_u(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int o = m.o, v = m.v;
    GRID_LOOP(e, (long long)o * v * o * v) {
        int b = (int)(e % v);
        long long r = e / v;
        int j = (int)(r % o); r /= o;
        int a = (int)(r % v);
        int i = (int)(r / v);
        m.u[e] = 2.0 * m.t2[e] - m.t2[(((long long)i * v + b) * o + j) * v + a];
    }
}

// Ts[i][mu][j][nu] *= G[mu][nu]
__global__ void k_gamma_scale(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int n = m.N, o = m.o;
    GRID_LOOP(e, (long long)o * n * o * n) {
        int nu = (int)(e % n);
        int mu = (int)((e / ((long long)n * o)) % n);
        m.Ts[e] *= m.G[mu * n + nu];
    }
}

// r1[i][a] = Fd[o+a][i];  Fvv2 = Fd_vv;  Foo2 = Fd_oo
__global__ void k_fock_blocks(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int n = m.N, o = m.o, v = m.v;
    GRID_LOOP(e, (long long)o * v + v * v + o * o) {
        if (e < o * v) {
            int i = (int)(e / v), a = (int)(e % v);
            m.r1[e] = m.Fd[(o + a) * n + i];
        } else if (e < o * v + v * v) {
            int f = (int)(e - o * v), b = f / v, c = f % v;
            m.Fvv2[f] = m.Fd[(o + b) * n + o + c];
        } else {
            int f = (int)(e - o * v - v * v), k = f / o, j = f % o;
            m.Foo2[f] = m.Fd[k * n + j];
        }
    }
}

// X2[i][a][j][b] = 0.5 Cp[i][a][j][b] + Cp[j][a][i][b]
__global__ void k_c_combine(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int o = m.o, v = m.v;
    GRID_LOOP(e, (long long)o * v * o * v) {
        int b = (int)(e % v);
        long long r = e / v;
        int j = (int)(r % o); r /= o;
        int a = (int)(r % v);
        int i = (int)(r / v);
        m.X2[e] = 0.5 * m.Cp[e] + m.Cp[(((long long)j * v + a) * o + i) * v + b];
    }
}

// r2 += X2 + X2^T (pair transpose)
__global__ void k_assemble(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const long long ov = (long long)m.o * m.v;
    GRID_LOOP(e, ov * ov) {
        long long p = e / ov, q = e % ov;
        m.r2[e] += m.X2[e] + m.X2[q * ov + p];
    }
}

// ---------------------------------------------------------------- step
// d1 = r1, d2 = 2 r2(ijab) - r2(ijba); t1 += s1 d1/D1 and, by the projection
// type of stepCC (mod_cc.f90:1007-1008),
//   "2-1" (proj 2): t2 += s2 (2 d2(ijab) + d2(ijba))/D2 = 3 s2 r2/D2,
//   "1"   (proj 1): t2 += s2 d2(ijab)/D2.
// Writes the new amplitudes and the DIIS error vector (d1, 3 r2 or d2, as
// pushCCVectors :1417-1420) into the history slot `slot`, and per-block
// maxima of |d1|, |d2| into part.
__global__ void k_step(const CCMol *mols, const DiisMol *diis, const int *active, double s1, double s2,
                       int use_diis, int proj, double *part, int nblk)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const DiisMol &h = diis[blockIdx.y];
    const int o = m.o, v = m.v;
    const long long ov = (long long)o * v, L2 = ov * ov;
    const int slot = h.count[0] % h.nd;
    double *Ht = use_diis ? h.Ht + (long long)slot * h.L : nullptr;
    double *He = use_diis ? h.He + (long long)slot * h.L : nullptr;
    double mx1 = 0.0, mx2 = 0.0;
    GRID_LOOP(e, ov + L2) {
        if (e < ov) {
            double d = m.r1[e];
            mx1 = fmax(mx1, fabs(d));
            double t = m.t1[e] + s1 * d / m.D1[e];
            m.t1[e] = t;
            if (Ht) { Ht[e] = t; He[e] = d; }
        } else {
            long long f = e - ov;
            int b = (int)(f % v);
            long long r = f / v;
            int j = (int)(r % o); r /= o;
            int a = (int)(r % v);
            int i = (int)(r / v);
            // as the reference, each pair (ia),(jb) takes the value computed for
            // (ia) <= (jb), so the amplitudes stay exactly pair-symmetric
            const long long p1 = (long long)i * v + a, q1 = (long long)j * v + b;
            const long long p2 = (long long)i * v + b, q2 = (long long)j * v + a;
            double w = m.r2[min(p1, q1) * ov + max(p1, q1)];
            double d2 = 2.0 * w - m.r2[min(p2, q2) * ov + max(p2, q2)];
            mx2 = fmax(mx2, fabs(d2));
            const double g = proj == 1 ? d2 : 3.0 * w;
            double t = m.t2[f] + s2 * g / m.D2[f];
            m.t2[f] = t;
            if (Ht) { Ht[e] = t; He[e] = g; }
        }
    }
    double r1 = block_red(mx1, true);
    double r2 = block_red(mx2, true);
    if (threadIdx.x == 0) {
        part[((long long)blockIdx.y * nblk + blockIdx.x) * 2 + 0] = r1;
        part[((long long)blockIdx.y * nblk + blockIdx.x) * 2 + 1] = r2;
    }
}

__global__ void k_step_finish(const CCMol *mols, const int *active, const double *part, int nblk)
{
    const int mol = blockIdx.x;
    if (active && !active[mol]) return;
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
        a = fmax(a, part[((long long)mol * nblk + k) * 2 + 0]);
        b = fmax(b, part[((long long)mol * nblk + k) * 2 + 1]);
    }
    a = warp_max(a); b = warp_max(b);
    if (threadIdx.x == 0) { mols[mol].res[0] = a; mols[mol].res[1] = b; }
}

// ---------------------------------------------------------------- DIIS
// gate[mol]: the DIIS step runs while max(|d1|,|d2|) >= gate[mol]. The
// reference stops mixing once the residual is below the convergence target
// (there the iteration ends); FP64 iterations use that target, tensor-core
// iterations (which hand over rather than converge) their hand-over target.
// Weighted dots of the newest error vector with every stored one. The doubles
// part is a symmetric pair matrix; the reference's vectors hold only the pairs
// (ia) <= (jb), so off-diagonal products count 1/2 and diagonal ones 1.
__global__ void k_diis_dots(const CCMol *mols, const DiisMol *diis, const int *active, const double *gate,
                            double *part, int nblk)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const DiisMol &h = diis[blockIdx.y];
    if (!(fmax(m.res[0], m.res[1]) >= gate[blockIdx.y])) return;      // converged: the reference skips DIIS
    const long long ov = (long long)m.o * m.v;
    const int cnt = h.count[0] + 1, n = cnt < h.nd ? cnt : h.nd;
    const int k = blockIdx.z;                             // stored vector of this block
    if (k >= n) return;
    const int slot = h.count[0] % h.nd;
    const double *en = h.He + (long long)slot * h.L;
    const double *ek = h.He + (long long)k * h.L;
    double acc = 0.0;
    GRID_LOOP(e, h.L) {
        double w = 1.0;
        if (e >= ov) {
            long long f = e - ov, p = f / ov, q = f % ov;
            w = (p == q) ? 1.0 : 0.5;
        }
        acc += w * en[e] * ek[e];
    }
    double r = block_red(acc, false);
    if (threadIdx.x == 0) part[((long long)blockIdx.y * nblk + blockIdx.x) * HX_MAX_DIIS + k] = r;
}

// Ordered sum of the partial dots into the Gram matrix (slot indexing), then
// the bordered DIIS system solved by Gaussian elimination with partial
// pivoting (one thread per molecule). Coefficients go to h.coef[slot].
__global__ void k_diis_solve(const CCMol *mols, const DiisMol *diis, const int *active, const double *gate,
                             const double *part, int nblk)
{
    const int mol = blockIdx.x;
    if (active && !active[mol]) return;
    const CCMol &m = mols[mol];
    const DiisMol &h = diis[mol];
    if (!(fmax(m.res[0], m.res[1]) >= gate[mol])) return;
    const int cnt = h.count[0] + 1, n = cnt < h.nd ? cnt : h.nd;
    const int slot = h.count[0] % h.nd;
    __shared__ double g[HX_MAX_DIIS];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += part[((long long)mol * nblk + b) * HX_MAX_DIIS + k];
        g[k] = s;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int k = 0; k < n; ++k) {
        h.gram[slot * h.nd + k] = g[k];
        h.gram[k * h.nd + slot] = g[k];
    }
    h.count[0] = cnt;
    if (n == 1) { h.coef[HX_MAX_DIIS] = 0.0; return; }     // newCCVectors(1) returns early
    const int nb = n + 1;
    double A[(HX_MAX_DIIS + 1) * (HX_MAX_DIIS + 1)], x[HX_MAX_DIIS + 1];
    for (int p = 0; p < nb; ++p) {
        for (int q = 0; q < nb; ++q) {
            double val;
            if (p == n && q == n) val = 0.0;
            else if (p == n || q == n) val = 1.0;
            else val = h.gram[p * h.nd + q];
            A[p * nb + q] = val;
        }
        x[p] = (p == n) ? 1.0 : 0.0;
    }
    for (int k = 0; k < nb; ++k) {
        int piv = k;
        for (int r = k + 1; r < nb; ++r)
            if (fabs(A[r * nb + k]) > fabs(A[piv * nb + k])) piv = r;
        if (piv != k) {
            for (int c = 0; c < nb; ++c) { double t = A[k * nb + c]; A[k * nb + c] = A[piv * nb + c]; A[piv * nb + c] = t; }
            double t = x[k]; x[k] = x[piv]; x[piv] = t;
        }
        for (int r = k + 1; r < nb; ++r) {
            double f = A[r * nb + k] / A[k * nb + k];
            for (int c = k; c < nb; ++c) A[r * nb + c] -= f * A[k * nb + c];
            x[r] -= f * x[k];
        }
    }
    for (int k = nb - 1; k >= 0; --k) {
        double s = x[k];
        for (int c = k + 1; c < nb; ++c) s -= A[k * nb + c] * x[c];
        x[k] = s / A[k * nb + k];
    }
    for (int k = 0; k < n; ++k) {
        if (!isfinite(x[k])) { h.coef[HX_MAX_DIIS] = 0.0; return; }   // singular subspace: no mixing
        h.coef[k] = x[k];
    }
    h.coef[HX_MAX_DIIS] = (double)n;     // number of vectors to mix
}

// t = sum_k c_k Ht[k]
__global__ void k_diis_extrapolate(const CCMol *mols, const DiisMol *diis, const int *active, const double *gate)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const DiisMol &h = diis[blockIdx.y];
    if (!(fmax(m.res[0], m.res[1]) >= gate[blockIdx.y])) return;
    const int n = (int)h.coef[HX_MAX_DIIS];
    if (n < 2) return;
    const long long ov = (long long)m.o * m.v;
    GRID_LOOP(e, h.L) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += h.coef[k] * h.Ht[(long long)k * h.L + e];
        if (e < ov) m.t1[e] = s; else m.t2[e - ov] = s;
    }
}

// ---------------------------------------------------------------- energy
// E = 2 sum F_ia t_ia + sum_(ia),(jb) L(ia,jb) (t2 + t1 t1)   (energyCC r-ccsd)
__global__ void k_energy(const CCMol *mols, const int *active, double *part, int nblk)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int o = m.o, v = m.v, n = m.N;
    const long long ov = (long long)o * v;
    double s1 = 0.0, s2 = 0.0;
    GRID_LOOP(e, ov + ov * ov) {
        if (e < ov) {
            int i = (int)(e / v), a = (int)(e % v);
            s1 += m.Fmo[i * n + o + a] * m.t1[e];
        } else {
            long long f = e - ov, p = f / ov, q = f % ov;
            s2 += m.Lov[f] * (m.t2[f] + m.t1[p] * m.t1[q]);
        }
    }
    double r1 = block_red(s1, false);
    double r2 = block_red(s2, false);
    if (threadIdx.x == 0) {
        part[((long long)blockIdx.y * nblk + blockIdx.x) * 2 + 0] = r1;
        part[((long long)blockIdx.y * nblk + blockIdx.x) * 2 + 1] = r2;
    }
}

__global__ void k_energy_finish(const CCMol *mols, const int *active, const double *part, int nblk)
{
    const int mol = blockIdx.x;
    if (active && !active[mol]) return;
    if (threadIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nblk; ++k) {
        a += part[((long long)mol * nblk + k) * 2 + 0];
        b += part[((long long)mol * nblk + k) * 2 + 1];
    }
    const CCMol &m = mols[mol];
    m.res[2] = 2.0 * a + b + m.eref;
    m.res[3] = m.eref;
    m.res[4] = 2.0 * a;
    m.res[5] = b;
}

// ---------------------------------------------------------------- set-up
// Constants after SCF: denominators, ZDO vectors of the undressed ov space,
// and the reference guess (guessCC r-ccsd, mod_cc.f90:634-650) when asked.
__global__ void k_setup(const CCMol *mols, const int *active)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int n = m.N, o = m.o, v = m.v;
    const long long ov = (long long)o * v;
    GRID_LOOP(e, ov + ov * ov + (long long)n * ov) {
        if (e < ov) {
            int i = (int)(e / v), a = (int)(e % v);
            m.D1[e] = m.Fmo[i * n + i] - m.Fmo[(o + a) * n + o + a];
        } else if (e < ov + ov * ov) {
            long long f = e - ov;
            int b = (int)(f % v);
            long long r = f / v;
            int j = (int)(r % o); r /= o;
            int a = (int)(r % v);
            int i = (int)(r / v);
            // grouped so that (ia),(jb) and (jb),(ia) round identically
            m.D2[f] = (m.Fmo[i * n + i] + m.Fmo[j * n + j]) - (m.Fmo[(o + a) * n + o + a] + m.Fmo[(o + b) * n + o + b]);
        } else {
            long long f = e - ov - ov * ov;
            int mu = (int)(f / ov), r = (int)(f % ov), k = r / v, c = r % v;
            m.Bov0[f] = m.Cmo[mu * n + k] * m.Cmo[mu * n + o + c];
        }
    }
}

// Lov = 2 gov - gov(ab swapped); t1, t2 = reference guess (when guess != 0)
__global__ void k_setup2(const CCMol *mols, const int *active, int guess)
{
    if (skip(active)) return;
    const CCMol &m = mols[blockIdx.y];
    const int n = m.N, o = m.o, v = m.v;
    const long long ov = (long long)o * v;
    GRID_LOOP(e, ov * ov) {
        int b = (int)(e % v);
        long long r = e / v;
        int j = (int)(r % o); r /= o;
        int a = (int)(r % v);
        int i = (int)(r / v);
        // canonical (upper-triangle) values: the guess and L are exactly pair-symmetric
        const long long p1 = (long long)i * v + a, q1 = (long long)j * v + b;
        const long long p2 = (long long)i * v + b, q2 = (long long)j * v + a;
        double g = m.gov[min(p1, q1) * ov + max(p1, q1)];
        double gx = m.gov[min(p2, q2) * ov + max(p2, q2)];
        double L = 2.0 * g - gx;
        m.Lov[e] = L;
        if (guess) m.t2[e] = L / m.D2[e];     // R(i,a,j,b) / (F_ii+F_jj-F_aa-F_bb)
        if (guess && e < ov) {
            int ii = (int)(e / v), aa = (int)(e % v);
            m.t1[e] = m.Fmo[ii * n + o + aa] / m.D1[e];
        }
    }
}
}  // namespace

// ---------------------------------------------------------------- launchers
static inline dim3 grid_for(long long work, int nmol, int cap = 4096)
{
    long long b = (work + NT - 1) / NT;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return dim3((unsigned)b, (unsigned)nmol);
}

#define LAUNCH_EW(kern, work, ...)                                                   \
    do {                                                                             \
        kern<<<grid_for(work, nmol), NT, 0, s>>>(__VA_ARGS__);                       \
        hx_count_launches(1);                                                        \
        cudaError_t e_ = cudaGetLastError();                                         \
        if (e_ != cudaSuccess) return e_;                                            \
    } while (0)

cudaError_t hx_ew_dress_init(const CCMol *m, const int *act, int nmol, long long maxw, cudaStream_t s)
{ LAUNCH_EW(k_dress_init, maxw, m, act); return cudaSuccess; }
cudaError_t hx_ew_dress_fock(const CCMol *m, const int *act, int nmol, long long maxw, cudaStream_t s)
{ LAUNCH_EW(k_dress_fock, maxw, m, act); return cudaSuccess; }
cudaError_t hx_ew_zdo_products(const CCMol *m, const int *act, int nmol, long long maxw, cudaStream_t s)
{ LAUNCH_EW(k_zdo_products, maxw, m, act); return cudaSuccess; }
cudaError_t hx_ew_make_u(const CCMol *m, const int *act, int nmol, long long maxw, cudaStream_t s)
{ LAUNCH_EW(k_make_u, maxw, m, act); return cudaSuccess; }
cudaError_t hx_ew_gamma_scale(const CCMol *m, const int *act, int nmol, long long maxw, cudaStream_t s)
{ LAUNCH_EW(k_gamma_scale, maxw, m, act); return cudaSuccess; }
cudaError_t hx_ew_fock_blocks(const CCMol *m, const int *act, int nmol, long long maxw, cudaStream_t s)
{ LAUNCH_EW(k_fock_blocks, maxw, m, act); return cudaSuccess; }
cudaError_t hx_ew_c_combine(const CCMol *m, const int *act, int nmol, long long maxw, cudaStream_t s)
{ LAUNCH_EW(k_c_combine, maxw, m, act); return cudaSuccess; }
cudaError_t hx_ew_assemble(const CCMol *m, const int *act, int nmol, long long maxw, cudaStream_t s)
{ LAUNCH_EW(k_assemble, maxw, m, act); return cudaSuccess; }
cudaError_t hx_ew_setup(const CCMol *m, const int *act, int nmol, long long maxw, int guess, cudaStream_t s)
{
    LAUNCH_EW(k_setup, maxw, m, act);
    return cudaSuccess;
}
cudaError_t hx_ew_setup2(const CCMol *m, const int *act, int nmol, long long maxw, int guess, cudaStream_t s)
{
    LAUNCH_EW(k_setup2, maxw, m, act, guess);
    return cudaSuccess;
}

cudaError_t hx_step(const CCMol *m, const DiisMol *h, const int *act, int nmol, double s1, double s2,
                    int use_diis, int proj, double *part, int nblk, cudaStream_t s)
{
    k_step<<<dim3(nblk, nmol), NT, 0, s>>>(m, h, act, s1, s2, use_diis, proj, part, nblk);
    hx_count_launches(2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_step_finish<<<nmol, 32, 0, s>>>(m, act, part, nblk);
    return cudaGetLastError();
}

cudaError_t hx_diis(const CCMol *m, const DiisMol *h, const int *act, int nmol, const double *gate, double *part,
                    int nblk, int nd_max, cudaStream_t s)
{
    k_diis_dots<<<dim3(nblk, nmol, nd_max), NT, 0, s>>>(m, h, act, gate, part, nblk);
    hx_count_launches(3);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_diis_solve<<<nmol, 32, 0, s>>>(m, h, act, gate, part, nblk);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_diis_extrapolate<<<dim3(nblk, nmol), NT, 0, s>>>(m, h, act, gate);
    return cudaGetLastError();
}

cudaError_t hx_energy(const CCMol *m, const int *act, int nmol, double *part, int nblk, cudaStream_t s)
{
    k_energy<<<dim3(nblk, nmol), NT, 0, s>>>(m, act, part, nblk);
    hx_count_launches(2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_energy_finish<<<nmol, 32, 0, s>>>(m, act, part, nblk);
    return cudaGetLastError();
}
