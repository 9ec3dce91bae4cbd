// Elementwise, reduction and DIIS kernels of the CCSD iteration (FP64, HBM bound).
//
// All kernels are grouped over the molecules of a batch with a balanced
// schedule (HxSched, hx_plan.h): every molecule owns a run of blocks in
// proportion to its work, a block finds its molecule by binary search over
// the prefix sums, and blocks of molecules whose `active` flag is 0 return at
// once. Reductions are two-pass (fixed per-block partials, then an ordered
// sum per molecule), so repeated runs are bitwise identical.
//
// The amplitude tail of an iteration (stepCC, pushCCVectors, diisDotProduct,
// newCCVectors and energyCC; mod_cc.f90:987-1017, 1390-1423, 1514-1555,
// 2133-2193, 1916-1952) works on "pair units": v x v blocks [a][b] of the
// pair matrix for occupied pairs (i, j), staged in shared memory so that the
// (a, b) transposes the equations need are read and written coalesced.
//   k_step_push   residual assembly (r2 + X2 + X2 pair-transposed), the
//                 Jacobi step, the push into the DIIS ring and the dots of
//                 the new error vector with every stored one, per unit;
//   k_diis_solve  per molecule: maxima, Gram row, bordered solve;
//   k_extrapolate t = sum c_k t_k written to both halves of t2, and the
//                 energy partials of the result.
// Only the canonical blocks i <= j are stepped and stored, as the reference
// stores only the pairs (ia) <= (jb).
#include "hx_common.cuh"
#include "hx_plan.h"
#include "hx_kernels.h"

namespace {
constexpr int NT = 256;

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
// block-wide reduction (sum or max) of blockDim.x == NT threads; the result is
// valid in thread 0 and the shared scratch may be reused after the call
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
    return v;
}

// molecule of block b: the last m with start[m] <= b
__device__ __forceinline__ int sched_mol(const int *__restrict__ start, int nmol, int b)
{
    int lo = 0, hi = nmol - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Element-wise kernels: block b of molecule mol covers HX_EW_CHUNK elements.
#define EW_PROLOGUE                                                                      \
    const int mol_ = sched_mol(start, nmol, blockIdx.x);                                 \
    if (active && !active[mol_]) return;                                                 \
    const CCMol &m = mols[mol_];                                                         \
    const long long base_ = (long long)(blockIdx.x - start[mol_]) * HX_EW_CHUNK;
#define EW_LOOP(e, n)                                                                    \
    for (long long e = base_ + threadIdx.x, end_ = min(base_ + HX_EW_CHUNK, (long long)(n)); e < end_; e += NT)
#define EW_ARGS const CCMol *__restrict__ mols, const int *__restrict__ active, const int *__restrict__ start, int nmol

// ---------------------------------------------------------------- dressing
// X = [Co | Cv], Y = [Co | Cv]; the t1 corrections are added by GEMMs.
__global__ void k_dress_init(EW_ARGS)
{
    EW_PROLOGUE
    EW_LOOP(e, (long long)m.N * m.N) { m.X[e] = m.Cmo[e]; m.Y[e] = m.Cmo[e]; }
}

// H2 = h - G o Pm + 2 diag(G diag Pm), Pm = Yo Xo^T (dressed half density)
__global__ void k_dress_fock(EW_ARGS)
{
    EW_PROLOGUE
    const int n = m.N;
    EW_LOOP(e, (long long)n * n) {
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
__global__ void k_zdo_products(EW_ARGS)
{
    EW_PROLOGUE
    const int n = m.N, o = m.o, v = m.v;
    const long long nia = (long long)n * o * v, noo = (long long)n * o * o, nvv = (long long)n * v * v;
    EW_LOOP(e, nia + noo + nvv) {
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

// Ts[i][mu][j][nu] *= G[mu][nu]  (a molecule's o N o N < 2^32 elements: 32-bit index arithmetic)
__global__ void k_gamma_scale(EW_ARGS)
{
    EW_PROLOGUE
    const unsigned n = (unsigned)m.N, no = n * (unsigned)m.o;
    double *__restrict__ Ts = m.Ts;
    const double *__restrict__ G = m.G;
    EW_LOOP(e, (long long)no * no) {
        const unsigned x = (unsigned)e;
        const unsigned nu = x % n, mu = (x / no) % n;
        Ts[e] *= G[mu * n + nu];
    }
}

// r1[i][a] = Fd[o+a][i];  Fvv2 = Fd_vv;  Foo2 = Fd_oo
__global__ void k_fock_blocks(EW_ARGS)
{
    EW_PROLOGUE
    const int n = m.N, o = m.o, v = m.v;
    EW_LOOP(e, (long long)o * v + v * v + o * o) {
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

// X2[i][a][j][b] = 0.5 Cp[i][a][j][b] + Cp[j][a][i][b]  (consecutive b read consecutively)
__global__ void k_c_combine(EW_ARGS)
{
    EW_PROLOGUE
    const unsigned o = (unsigned)m.o, v = (unsigned)m.v;
    const double *__restrict__ Cp = m.Cp;
    double *__restrict__ X2 = m.X2;
    EW_LOOP(e, (long long)o * v * o * v) {
        const unsigned x = (unsigned)e;                  // o^2 v^2 < 2^32
        const unsigned b = x % v, r = x / v, j = r % o, r2 = r / o, a = r2 % v, i = r2 / v;
        X2[e] = 0.5 * Cp[e] + Cp[((j * v + a) * o + i) * v + b];
    }
}

// ---------------------------------------------------------------- pair units
// Units of one molecule: unit 0 is the singles; unit u >= 1 holds the v x v
// blocks [(u-1) g, min(u g, nb)) of the occupied pairs (i, j), in row-major
// order of the upper triangle i <= j (SK_UP) or of the whole o x o grid
// (SK_FULL), g = hx_unit_blocks(v). A unit's blocks sit in shared memory as
// [block][a][b] with rows padded to v + 1 (transposed reads spread over banks).
struct Unit {
    int mol, u, k0, nb;   // molecule, unit, first block, blocks in this unit
};

// (i, j) of block k of the upper triangle (row i starts at i o - i (i - 1) / 2)
__device__ __forceinline__ void up_block(int k, int o, int &i, int &j)
{
    const double s = 2.0 * o + 1.0;
    int r = (int)((s - sqrt(s * s - 8.0 * k)) * 0.5);
    r = r < 0 ? 0 : (r > o - 1 ? o - 1 : r);
    while (r > 0 && r * o - r * (r - 1) / 2 > k) --r;
    while (r + 1 < o && (r + 1) * o - (r + 1) * r / 2 <= k) ++r;
    i = r;
    j = r + (k - (r * o - r * (r - 1) / 2));
}

// This block's unit, and the (i, j) of its pair blocks in bi/bj (shared).
__device__ __forceinline__ Unit unit_of(const CCMol *mols, const int *start, int nmol, bool upper, int *bi, int *bj)
{
    Unit w;
    w.mol = sched_mol(start, nmol, blockIdx.x);
    w.u = blockIdx.x - start[w.mol];
    const CCMol &m = mols[w.mol];
    const int g = hx_unit_blocks(m.v);
    const int nbt = upper ? m.o * (m.o + 1) / 2 : m.o * m.o;
    w.k0 = w.u > 0 ? (w.u - 1) * g : 0;
    w.nb = w.u > 0 ? min(g, nbt - w.k0) : 0;
    for (int lb = threadIdx.x; lb < w.nb; lb += blockDim.x) {
        int i, j;
        if (upper) up_block(w.k0 + lb, m.o, i, j);
        else { i = (w.k0 + lb) / m.o; j = (w.k0 + lb) % m.o; }
        bi[lb] = i;
        bj[lb] = j;
    }
    __syncthreads();
    return w;
}

__device__ __forceinline__ long long pair_off(int i, int a, int j, int b, int o, int v)
{
    return (((long long)i * v + a) * o + j) * v + b;
}

// Tile loops of a unit: warp w walks the rows (block lb, row a) of the unit's
// tile, its lanes the columns b, so global reads and writes run along b (one
// division per row, none per element); shared-memory index of (lb, a, b) is
// (lb v + a)(v + 1) + b.
#define ROW_LOOP(nrows) for (int row_ = threadIdx.x >> 5; row_ < (nrows); row_ += NT / 32)
#define COL_LOOP(b, v) for (int b = threadIdx.x & 31; b < (v); b += 32)

// K sums over the block at once (two barriers); valid in thread 0
template <int K>
__device__ __forceinline__ void block_sum_n(double (&x)[K])
{
    __shared__ double sh[K][NT / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) x[k] = warp_sum(x[k]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) sh[k][w] = x[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        x[k] = (threadIdx.x < NT / 32) ? sh[k][threadIdx.x] : 0.0;
        if (w == 0) x[k] = warp_sum(x[k]);
    }
}

// u[i][a][j][b] = 2 t[i][a][j][b] - t[i][b][j][a]  (SK_FULL units)
__global__ void __launch_bounds__(NT) k_make_u(const CCMol *__restrict__ mols, const int *__restrict__ active,
                                               const int *__restrict__ start, int nmol)
{
    extern __shared__ double sm[];
    __shared__ int bi[64], bj[64];
    const Unit w = unit_of(mols, start, nmol, false, bi, bj);
    if ((active && !active[w.mol]) || w.u == 0) return;
    const CCMol &m = mols[w.mol];
    const int o = m.o, v = m.v, nrows = w.nb * v;
    const double *__restrict__ t2 = m.t2;
    double *__restrict__ u = m.u;
#pragma unroll 4
    ROW_LOOP(nrows) {
        const int lb = row_ / v, a = row_ - lb * v;
        const double *src = t2 + pair_off(bi[lb], a, bj[lb], 0, o, v);
        double *srow = sm + (lb * v + a) * (v + 1);
        COL_LOOP(b, v) srow[b] = src[b];
    }
    __syncthreads();
#pragma unroll 4
    ROW_LOOP(nrows) {
        const int lb = row_ / v, a = row_ - lb * v;
        double *dst = u + pair_off(bi[lb], a, bj[lb], 0, o, v);
        const double *srow = sm + (lb * v + a) * (v + 1);
        COL_LOOP(b, v) dst[b] = 2.0 * srow[b] - sm[(lb * v + b) * (v + 1) + a];
    }
}

// Residual, Jacobi step and DIIS push of one unit (SK_UP units).
//   singles: d1 = r1; t1 += s1 d1 / D1.
//   doubles of a block (i, j), i <= j: w = Omega2(ia, jb) assembled as
//     r2 + X2 + X2 pair-transposed (the E and C/D terms), d2 = 2 w(ab) - w(ba)
//     (= w on a diagonal block, whose canonical element is the same for both);
//     g = 3 w ("2-1") or d2 ("1"); t2 += s2 g / D2 with D2 = (F_ii + F_jj) -
//     (F_aa + F_bb) (the grouping the set-up uses, so (ia,jb) and (jb,ia)
//     round alike).
// push = 1: (t, g) go into the ring slot count % nd and part gets the dots of
// g with every stored error vector. The error vector keeps the pair (ia, ib)
// of a diagonal block once (a <= b; the mirror element is stored as 0), so a
// plain dot is the reference's packed dot over (ia) <= (jb); t2 itself is
// written by k_amplitudes_energy. push = 0 (no DIIS): t1 and both halves of t2 are
// written here. part[0], part[1] = max|d1|, max|d2|.
__global__ void __launch_bounds__(NT) k_step_push(const CCMol *__restrict__ mols, const DiisMol *__restrict__ diis,
                                                  const int *__restrict__ active, const int *__restrict__ start,
                                                  int nmol, double s1, double s2, int proj, int push,
                                                  double *__restrict__ part)
{
    extern __shared__ double sm[];
    __shared__ int bi[64], bj[64];
    const Unit w = unit_of(mols, start, nmol, true, bi, bj);
    if (active && !active[w.mol]) return;
    const CCMol &m = mols[w.mol];
    const DiisMol &h = diis[w.mol];
    const int o = m.o, v = m.v, n = m.N, ov = o * v;
    double *P = part + (long long)blockIdx.x * HX_PART_STRIDE;
    const int cnt = push ? h.count[0] : 0;
    const int slot = push ? cnt % h.nd : 0, nvec = push ? min(cnt + 1, h.nd) : 0;
    const double *__restrict__ Fmo = m.Fmo;
    double *__restrict__ t2 = m.t2;
    const double *__restrict__ X2 = m.X2;
    double *S = sm;                              // the assembled residual of the unit's blocks
    double mx = 0.0;
    long long hoff;
    const int nrows = w.nb * v;
    if (w.u == 0) {
        hoff = 0;
        for (int e = threadIdx.x; e < ov; e += NT) {
            const double d = m.r1[e];
            mx = fmax(mx, fabs(d));
            const double t = m.t1[e] + s1 * d / m.D1[e];
            if (push) { h.Ht[(long long)slot * h.L + e] = t; h.He[(long long)slot * h.L + e] = d; }
            else m.t1[e] = t;
        }
    } else {
        hoff = ov + (long long)w.k0 * v * v;
        // S = r2 + (X2 + X2[q][p]): element (a, b) of block (i, j) takes X2[j][b][i][a],
        // read along a (coalesced) and added at the transposed tile position
#pragma unroll 4
        ROW_LOOP(nrows) {
            const int lb = row_ / v, a = row_ - lb * v;
            const double *src = X2 + pair_off(bi[lb], a, bj[lb], 0, o, v);
            double *srow = S + (lb * v + a) * (v + 1);
            COL_LOOP(b, v) srow[b] = src[b];
        }
        __syncthreads();
#pragma unroll 4
        ROW_LOOP(nrows) {
            const int lb = row_ / v, x = row_ - lb * v;              // x plays b
            const double *src = X2 + pair_off(bj[lb], x, bi[lb], 0, o, v);
            COL_LOOP(y, v) S[(lb * v + y) * (v + 1) + x] += src[y];  // y plays a
        }
        __syncthreads();
#pragma unroll 4
        ROW_LOOP(nrows) {
            const int lb = row_ / v, a = row_ - lb * v;
            const double *src = m.r2 + pair_off(bi[lb], a, bj[lb], 0, o, v);
            double *srow = S + (lb * v + a) * (v + 1);
            COL_LOOP(b, v) srow[b] = src[b] + srow[b];
        }
        __syncthreads();
        ROW_LOOP(nrows) {
            const int lb = row_ / v, a = row_ - lb * v, i = bi[lb], j = bj[lb];
            const double fij = Fmo[i * n + i] + Fmo[j * n + j], faa = Fmo[(o + a) * n + o + a];
            const double *srow = S + (lb * v + a) * (v + 1);
            double *trow = t2 + pair_off(i, a, j, 0, o, v);
            const long long hrow = hoff + (long long)(lb * v + a) * v;
            COL_LOOP(b, v) {
                const double sab = srow[b], sba = S[(lb * v + b) * (v + 1) + a];
                double wv, d2;
                if (i < j) { wv = sab; d2 = 2.0 * sab - sba; }
                else { wv = a <= b ? sab : sba; d2 = wv; }
                mx = fmax(mx, fabs(d2));
                const double g = proj == 1 ? d2 : 3.0 * wv;
                const double D = fij - (faa + Fmo[(o + b) * n + o + b]);
                const double t = trow[b] + s2 * g / D;
                if (push) {
                    h.Ht[(long long)slot * h.L + hrow + b] = t;
                    // a diagonal block holds (ia, ib) and (ib, ia), the same pair: the
                    // error vector keeps it once (a <= b), so plain dots of stored error
                    // vectors are the reference's packed dots
                    h.He[(long long)slot * h.L + hrow + b] = (i == j && a > b) ? 0.0 : g;
                } else {
                    trow[b] = t;
                }
            }
        }
        __syncthreads();                         // (also makes the global writes above visible to the block)
        if (!push) {   // the mirror half: t2[j][b][i][a] = t2[i][a][j][b], a fastest (DIIS off only)
            ROW_LOOP(nrows) {
                const int lb = row_ / v, x = row_ - lb * v, i = bi[lb], j = bj[lb];   // x plays b
                if (i < j) {
                    double *dst = t2 + pair_off(j, x, i, 0, o, v);
                    COL_LOOP(y, v) dst[y] = t2[pair_off(i, y, j, x, o, v)];
                }
            }
        }
    }
    const double r = block_red(mx, true);
    if (threadIdx.x == 0) { P[0] = w.u == 0 ? r : 0.0; P[1] = w.u == 0 ? 0.0 : r; }
    // dots of the new error vector (just written, read back from L2) with every
    // stored one over the unit's contiguous stretch of the ring, eight stored
    // vectors per pass
    const int ne = w.u == 0 ? ov : w.nb * v * v;
    const double *En = h.He + (long long)slot * h.L + hoff;
    for (int k0 = 0; k0 < nvec; k0 += 8) {
        double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        const double *Ek[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) Ek[q] = h.He + (long long)(k0 + q < nvec ? k0 + q : slot) * h.L + hoff;
#pragma unroll 2
        for (int e = threadIdx.x; e < ne; e += NT) {
            const double g = En[e];
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[q] += g * Ek[q][e];
        }
        block_sum_n<8>(acc);
        if (threadIdx.x == 0)
            for (int q = 0; q < 8 && k0 + q < nvec; ++q) P[2 + k0 + q] = acc[q];
    }
}

// ---------------------------------------------------------------- DIIS
// One block per molecule. The maxima of the units give res[0], res[1] (the
// reference's accuracy(1..2), before the step). gate[mol]: the DIIS step runs
// while max(|d1|,|d2|) >= gate[mol]. The reference stops mixing once the
// residual is below the convergence target (there the iteration ends); FP64
// iterations use that target, tensor-core iterations (which hand over rather
// than converge) their hand-over target. When it runs, the units' dots
// summed in a fixed order (strided per thread, then a fixed tree) form the
// Gram row of the new slot and the bordered system is solved by Gaussian
// elimination with partial pivoting; coef[HX_MAX_DIIS] = vectors to mix (1:
// none, t = the newest) and coef[HX_MAX_DIIS + 1] = the newest slot.
__global__ void __launch_bounds__(NT) k_diis_solve(const CCMol *__restrict__ mols, const DiisMol *__restrict__ diis,
                                                   const int *__restrict__ active, const int *__restrict__ start,
                                                   const double *gate, const double *__restrict__ part, int push)
{
    const int mol = blockIdx.x;
    if (active && !active[mol]) return;
    const CCMol &m = mols[mol];
    const int u0 = start[mol], u1 = start[mol + 1];
    __shared__ double ab[2];
    double a = 0.0, b = 0.0;
    for (int u = u0 + threadIdx.x; u < u1; u += NT) {
        a = fmax(a, part[(long long)u * HX_PART_STRIDE + 0]);
        b = fmax(b, part[(long long)u * HX_PART_STRIDE + 1]);
    }
    a = block_red(a, true);
    b = block_red(b, true);
    if (threadIdx.x == 0) { m.res[0] = a; m.res[1] = b; ab[0] = a; ab[1] = b; }
    __syncthreads();
    a = ab[0];
    b = ab[1];
    if (!push) return;
    const DiisMol &h = diis[mol];
    const int cnt = h.count[0];
    const int slot = cnt % h.nd, n = cnt + 1 < h.nd ? cnt + 1 : h.nd;
    if (!(fmax(a, b) >= gate[mol])) {                  // converged: the reference skips DIIS
        if (threadIdx.x == 0) { h.coef[HX_MAX_DIIS] = 1.0; h.coef[HX_MAX_DIIS + 1] = slot; }
        return;
    }
    __shared__ double g[HX_MAX_DIIS];
    for (int k = 0; k < n; ++k) {
        double s = 0.0;
        for (int u = u0 + threadIdx.x; u < u1; u += NT) s += part[(long long)u * HX_PART_STRIDE + 2 + k];
        s = block_red(s, false);
        if (threadIdx.x == 0) g[k] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < n; ++k) {
            h.gram[slot * h.nd + k] = g[k];
            h.gram[k * h.nd + slot] = g[k];
        }
        h.count[0] = cnt + 1;
        h.coef[HX_MAX_DIIS + 1] = slot;
        h.coef[HX_MAX_DIIS] = 1.0;
    }
    if (n == 1) return;                                // newCCVectors(1) returns early
    // the bordered system [B 1; 1 0] c = e by Gaussian elimination with partial
    // pivoting in shared memory: pivot search and back substitution in one
    // thread, the row updates in parallel (each row's operations in the same
    // order as a serial elimination)
    constexpr int MB = HX_MAX_DIIS + 1;
    __shared__ double A[MB * MB], x[MB];
    __shared__ int piv_s;
    const int nb = n + 1;
    __syncthreads();
    for (int e = threadIdx.x; e < nb * nb; e += NT) {
        const int p = e / nb, q = e % nb;
        double val;
        if (p == n && q == n) val = 0.0;
        else if (p == n || q == n) val = 1.0;
        else val = h.gram[p * h.nd + q];
        A[p * nb + q] = val;
    }
    for (int p = threadIdx.x; p < nb; p += NT) x[p] = (p == n) ? 1.0 : 0.0;
    __syncthreads();
    for (int k = 0; k < nb; ++k) {
        if (threadIdx.x == 0) {
            int piv = k;
            for (int r = k + 1; r < nb; ++r)
                if (fabs(A[r * nb + k]) > fabs(A[piv * nb + k])) piv = r;
            piv_s = piv;
        }
        __syncthreads();
        const int piv = piv_s;
        if (piv != k) {
            for (int c = threadIdx.x; c < nb; c += NT) { double t = A[k * nb + c]; A[k * nb + c] = A[piv * nb + c]; A[piv * nb + c] = t; }
            if (threadIdx.x == 0) { double t = x[k]; x[k] = x[piv]; x[piv] = t; }
        }
        __syncthreads();
        for (int r = k + 1 + threadIdx.x; r < nb; r += NT) {
            const double f = A[r * nb + k] / A[k * nb + k];
            for (int c = k; c < nb; ++c) A[r * nb + c] -= f * A[k * nb + c];
            x[r] -= f * x[k];
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    for (int k = nb - 1; k >= 0; --k) {
        double s = x[k];
        for (int c = k + 1; c < nb; ++c) s -= A[k * nb + c] * x[c];
        x[k] = s / A[k * nb + k];
    }
    for (int k = 0; k < n; ++k)
        if (!isfinite(x[k])) return;                   // singular subspace: no mixing
    for (int k = 0; k < n; ++k) h.coef[k] = x[k];
    h.coef[HX_MAX_DIIS] = (double)n;
}

// ---------------------------------------------------------------- amplitudes and energy
// energyCC r-ccsd of the unit: part[0] = sum F_ia t_ia (singles unit),
// part[1] = the unit's share of sum L (t2 + t1 t1), where element (a, b) of
// block (i, j), i <= j, counts twice when i < j (it and its mirror) and once
// on a diagonal block. With DIIS (from != 0) the amplitudes come from the
// ring -- the newest vector, or sum_k c_k Ht[k] in slot order -- and are
// written to t1 and both halves of t2; without, they are read from t1, t2.
__global__ void __launch_bounds__(NT) k_amplitudes_energy(const CCMol *__restrict__ mols,
                                                          const DiisMol *__restrict__ diis,
                                                          const int *__restrict__ active,
                                                          const int *__restrict__ start, int nmol, int from,
                                                          double *__restrict__ part)
{
    extern __shared__ double sm[];
    __shared__ int bi[64], bj[64];
    __shared__ double cf[HX_MAX_DIIS];
    const Unit w = unit_of(mols, start, nmol, true, bi, bj);
    if (active && !active[w.mol]) return;
    const CCMol &m = mols[w.mol];
    const DiisMol &h = diis[w.mol];
    const int o = m.o, v = m.v, n = m.N, ov = o * v;
    const int nmix = from ? (int)h.coef[HX_MAX_DIIS] : 0, slot = from ? (int)h.coef[HX_MAX_DIIS + 1] : 0;
    for (int k = threadIdx.x; k < nmix; k += NT) cf[k] = h.coef[k];
    __syncthreads();
    const double *__restrict__ Ht = h.Ht;
    const long long L = h.L;
    auto combine = [&](long long e) {
        if (nmix <= 1) return Ht[(long long)slot * L + e];
        double s = 0.0;
#pragma unroll 4
        for (int k = 0; k < nmix; ++k) s += cf[k] * Ht[(long long)k * L + e];
        return s;
    };
    double *P = part + (long long)blockIdx.x * HX_PART_STRIDE;
    double acc = 0.0;
    double *__restrict__ t2 = m.t2;
    if (w.u == 0) {
        for (int e = threadIdx.x; e < ov; e += NT) {
            const double t = from ? combine(e) : m.t1[e];
            if (from) m.t1[e] = t;
            acc += m.Fmo[(e / v) * n + o + e % v] * t;
        }
    } else {
        // this unit's t1 rows i and j (from the ring: t1 is being written by unit 0)
        double *T1 = sm + hx_unit_tile(o, v);            // [block][2][v]
        for (int e = threadIdx.x; e < w.nb * 2 * v; e += NT) {
            const int lb = e / (2 * v), r = e % (2 * v), a = r % v, row = r < v ? bi[lb] : bj[lb];
            T1[e] = from ? combine((long long)row * v + a) : m.t1[row * v + a];
        }
        __syncthreads();
        const int nrows = w.nb * v;
        const long long hoff = ov + (long long)w.k0 * v * v;
#pragma unroll 2
        ROW_LOOP(nrows) {
            const int lb = row_ / v, a = row_ - lb * v, i = bi[lb], j = bj[lb];
            const long long f0 = pair_off(i, a, j, 0, o, v);
            double *trow = t2 + f0;
            const double *Lrow = m.Lov + f0;
            const double t1a = T1[lb * 2 * v + a];
            const long long hrow = hoff + (long long)(lb * v + a) * v;
            double *srow = sm + (lb * v + a) * (v + 1);
            COL_LOOP(b, v) {
                double t;
                if (from) {
                    t = combine(hrow + b);
                    trow[b] = t;
                    srow[b] = t;
                } else {
                    t = trow[b];
                }
                const double s = Lrow[b] * (t + t1a * T1[lb * 2 * v + v + b]);
                acc += i < j ? 2.0 * s : s;
            }
        }
        if (from) {
            __syncthreads();
            ROW_LOOP(nrows) {
                const int lb = row_ / v, x = row_ - lb * v, i = bi[lb], j = bj[lb];   // x plays b
                if (i < j) {
                    double *dst = t2 + pair_off(j, x, i, 0, o, v);
                    COL_LOOP(y, v) dst[y] = sm[(lb * v + y) * (v + 1) + x];
                }
            }
        }
    }
    const double r = block_red(acc, false);
    if (threadIdx.x == 0) { P[0] = w.u == 0 ? r : 0.0; P[1] = w.u == 0 ? 0.0 : r; }
}

// E = 2 sum F_ia t_ia + sum_(ia),(jb) L(ia,jb) (t2 + t1 t1)   (energyCC r-ccsd):
// the units' partials summed in a fixed order (strided per thread, fixed tree)
__global__ void __launch_bounds__(NT) k_energy_finish(const CCMol *__restrict__ mols, const int *__restrict__ active,
                                                      const int *__restrict__ start, const double *__restrict__ part)
{
    const int mol = blockIdx.x;
    if (active && !active[mol]) return;
    double x[2] = {0.0, 0.0};
    for (int u = start[mol] + threadIdx.x; u < start[mol + 1]; u += NT) {
        x[0] += part[(long long)u * HX_PART_STRIDE + 0];
        x[1] += part[(long long)u * HX_PART_STRIDE + 1];
    }
    block_sum_n<2>(x);
    if (threadIdx.x != 0) return;
    const CCMol &m = mols[mol];
    m.res[2] = 2.0 * x[0] + x[1] + m.eref;
    m.res[3] = m.eref;
    m.res[4] = 2.0 * x[0];
    m.res[5] = x[1];
}

// ---------------------------------------------------------------- set-up
// Constants after SCF: denominators, ZDO vectors of the undressed ov space,
// and the reference guess (guessCC r-ccsd, mod_cc.f90:634-650) when asked.
__global__ void k_setup(EW_ARGS)
{
    EW_PROLOGUE
    const int n = m.N, o = m.o, v = m.v;
    const long long ov = (long long)o * v;
    EW_LOOP(e, ov + ov * ov + (long long)n * ov) {
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
__global__ void k_setup2(EW_ARGS, int guess)
{
    EW_PROLOGUE
    const int n = m.N, o = m.o, v = m.v;
    const long long ov = (long long)o * v;
    EW_LOOP(e, ov * ov) {
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
#define LAUNCH_EW(kern, kind, ...)                                                                  \
    do {                                                                                            \
        if (S.blocks[kind] > 0)                                                                     \
            kern<<<(unsigned)S.blocks[kind], NT, 0, s>>>(m, act, S.start[kind], S.nmol, ##__VA_ARGS__); \
        hx_count_launches(1);                                                                       \
        cudaError_t e_ = cudaGetLastError();                                                        \
        if (e_ != cudaSuccess) return e_;                                                           \
    } while (0)

cudaError_t hx_ew_dress_init(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s)
{ LAUNCH_EW(k_dress_init, SK_NN); return cudaSuccess; }
cudaError_t hx_ew_dress_fock(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s)
{ LAUNCH_EW(k_dress_fock, SK_NN); return cudaSuccess; }
cudaError_t hx_ew_zdo_products(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s)
{ LAUNCH_EW(k_zdo_products, SK_ZDO); return cudaSuccess; }
cudaError_t hx_ew_gamma_scale(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s)
{ LAUNCH_EW(k_gamma_scale, SK_ONON); return cudaSuccess; }
cudaError_t hx_ew_fock_blocks(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s)
{ LAUNCH_EW(k_fock_blocks, SK_FOCK); return cudaSuccess; }
cudaError_t hx_ew_c_combine(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s)
{ LAUNCH_EW(k_c_combine, SK_PAIR); return cudaSuccess; }
cudaError_t hx_ew_setup(const CCMol *m, const int *act, const HxSched &S, cudaStream_t s)
{ LAUNCH_EW(k_setup, SK_SETUP); return cudaSuccess; }
cudaError_t hx_ew_setup2(const CCMol *m, const int *act, const HxSched &S, int guess, cudaStream_t s)
{ LAUNCH_EW(k_setup2, SK_PAIR, guess); return cudaSuccess; }

// dynamic shared memory of the pair-unit kernels (bytes): the largest over the batch
size_t hx_unit_smem(const int *o, const int *v, int nmol, int kernel)
{
    long long mx = 0;
    for (int k = 0; k < nmol; ++k) {
        const long long t = hx_unit_tile(o[k], v[k]);
        long long need = t;                                                 // k_make_u
        if (kernel == 1) need = t;                                          // k_step_push
        if (kernel == 2) need = t + 2LL * hx_unit_blocks(v[k]) * v[k];      // k_amplitudes_energy
        mx = need > mx ? need : mx;
    }
    return (size_t)mx * sizeof(double);
}

cudaError_t hx_unit_kernels_init(size_t smem_max)
{
    cudaError_t e = cudaSuccess;
    const int b = (int)smem_max;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_make_u, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_step_push, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_amplitudes_energy, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    return e;
}

cudaError_t hx_ew_make_u(const CCMol *m, const int *act, const HxSched &S, size_t smem, cudaStream_t s)
{
    k_make_u<<<(unsigned)S.blocks[SK_FULL], NT, smem, s>>>(m, act, S.start[SK_FULL], S.nmol);
    hx_count_launches(1);
    return cudaGetLastError();
}

// stepCC + pushCCVectors + diisDotProduct + newCCVectors + energyCC of every active molecule
cudaError_t hx_tail(const CCMol *m, const DiisMol *h, const int *act, const HxSched &S, const size_t smem[2],
                    double s1, double s2, int proj, int use_diis, const double *gate, double *part, cudaStream_t s)
{
    k_step_push<<<(unsigned)S.blocks[SK_UP], NT, smem[0], s>>>(m, h, act, S.start[SK_UP], S.nmol, s1, s2, proj,
                                                               use_diis, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_diis_solve<<<S.nmol, NT, 0, s>>>(m, h, act, S.start[SK_UP], gate, part, use_diis);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_amplitudes_energy<<<(unsigned)S.blocks[SK_UP], NT, smem[1], s>>>(m, h, act, S.start[SK_UP], S.nmol, use_diis,
                                                                       part);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_energy_finish<<<S.nmol, NT, 0, s>>>(m, act, S.start[SK_UP], part);
    hx_count_launches(4);
    return cudaGetLastError();
}

// energyCC of every (active) molecule from its current amplitudes
cudaError_t hx_energy(const CCMol *m, const DiisMol *h, const int *act, const HxSched &S, size_t smem, double *part,
                      cudaStream_t s)
{
    k_amplitudes_energy<<<(unsigned)S.blocks[SK_UP], NT, smem, s>>>(m, h, act, S.start[SK_UP], S.nmol, 0, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_energy_finish<<<S.nmol, NT, 0, s>>>(m, act, S.start[SK_UP], part);
    hx_count_launches(2);
    return cudaGetLastError();
}
